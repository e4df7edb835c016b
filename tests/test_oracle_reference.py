"""The CPU oracle against the reference's own generated code and FD checks.

The golden file holds outputs of the reference's symbolic derivative routines and
barrier functions (compiled from its sources by tests/golden/make_golden.py).
The finite-difference checks mirror the reference's derivTest_* and Check_*
routines (EDGE_EDGE_MOLLIFIER.h:384-580), using central differences.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_derivs.npz")
KIND = {"PE3D": 1, "PT": 2, "EE": 3, "EECN2": 4}


@pytest.mark.parametrize("name", ["PT", "EE", "PE3D", "EECN2"])
def test_derivatives_match_reference_generated_code(orc, name):
    z = np.load(GOLD)
    X, G, H = z["x_" + name], z["g_" + name], z["H_" + name]
    for x, g_ref, h_ref in zip(X, G, H):
        g, h = orc.d2_grad_hess(KIND[name], x)
        scale_g = np.abs(g_ref).max()
        scale_h = np.abs(h_ref).max()
        assert np.abs(g - g_ref).max() <= 1e-10 * scale_g
        # the generated Hessians are symmetric; storage order does not matter
        assert np.abs(h - h_ref).max() <= 1e-9 * scale_h


def test_barrier_matches_reference(orc):
    z = np.load(GOLD)
    for d, dhat, kappa, b, g, h in z["barrier"]:
        out = orc.barrier(d, dhat, kappa)
        for mine, ref in zip(out, (b, g, h)):
            assert abs(mine - ref) <= 1e-12 * max(abs(ref), 1e-300)


def test_elastic_barrier_is_offset_form_with_scaled_kappa(orc):
    # the reference's elastic-IPC barrier -kappa (s/shat - 1)^2 ln(s/shat) and its
    # derivatives equal the offset-IPC barrier with kappa / shat^2, the identity
    # the elastic-IPC path here is built on
    z = np.load(GOLD)
    for d, dhat, kappa, b, g, h in z["barrier_elastic"]:
        out = orc.barrier(d, dhat, kappa / (dhat * dhat))
        for mine, ref in zip(out, (b, g, h)):
            assert abs(mine - ref) <= 1e-12 * max(abs(ref), 1e-300), (d, dhat, mine, ref)


def test_strain_barrier_matches_reference(orc):
    # the strain-limiting barrier of one singular value against the reference's
    # f/g/h_sl_u (upper limit) and f/g/h_sl_l (lower limit) of INEXT.h, C2 form
    z = np.load(GOLD)
    rows = z["strain_barrier"]
    assert set(rows[:, 0]) == {0.0, 1.0}
    for _, sv, slim, shat, f, g, h in rows:
        out = orc.sl_barrier(sv, slim, shat)
        for mine, ref in zip(out, (f, g, h)):
            assert abs(mine - ref) <= 1e-13 * max(abs(ref), 1e-300), (sv, slim, shat, mine, ref)


def test_friction_mollifier_matches_reference(orc):
    # f0, f1 / |u| and the f2 term of the C1 friction mollifier against the
    # reference's FRICTION_UTILS.h on both sides of |u| = epsv h
    z = np.load(GOLD)
    rows = z["friction"]
    assert (rows[:, 0] < rows[:, 1] ** 2).any() and (rows[:, 0] >= rows[:, 1] ** 2).any()
    for x2, eh, f0, f1, f2 in rows:
        out = orc.friction_scalars(x2, eh)
        for mine, ref in zip(out, (f0, f1, f2)):
            assert abs(mine - ref) <= 1e-14 * abs(ref), (x2, eh, mine, ref)


def test_dihedral_angle_derivatives_match_reference(orc):
    # the reference's generated g_DA / H_DA differentiate the unsigned (acos)
    # angle; the bending energy uses the signed one, so they agree up to the sign
    # of the angle, (n2 x n1).(x1 - x2) with n1 = (x1-x0) x (x2-x0), n2 = (x2-x3) x (x1-x3)
    z = np.load(GOLD)
    signs = set()
    for x, g_ref, h_ref in zip(z["x_DA"], z["g_DA"], z["H_DA"]):
        v0, v1, v2, v3 = x[:3], x[3:6], x[6:9], x[9:]
        n1, n2 = np.cross(v1 - v0, v2 - v0), np.cross(v2 - v3, v1 - v3)
        sg = -1.0 if np.cross(n2, n1) @ (v1 - v2) < 0 else 1.0
        signs.add(sg)
        g, h = orc.dihedral_derivs(x)
        assert np.abs(g - sg * g_ref).max() <= 1e-11 * np.abs(g_ref).max()
        assert np.abs(h - sg * h_ref).max() <= 1e-9 * np.abs(h_ref).max()
    assert signs == {-1.0, 1.0}


def test_ee_mollifier_matches_reference(orc):
    # e(c) = (2 - c/eps) c/eps of c = |ea x eb|^2 below eps, with gradient and
    # Hessian by the chain rule, against the reference's EEM / g_EEM / H_EEM
    # composed with its g_EECN2 / H_EECN2
    z = np.load(GOLD)
    for x, eps, e_ref, g_ref, h_ref in zip(z["x_EEM"], z["eps_EEM"], z["e_EEM"], z["g_EEM"], z["H_EEM"]):
        e, g, h = orc.mollifier(x, eps)
        assert abs(e - e_ref) <= 1e-14 * abs(e_ref)
        assert np.abs(g - g_ref).max() <= 1e-10 * np.abs(g_ref).max()
        assert np.abs(h - h_ref).max() <= 1e-9 * np.abs(h_ref).max()


def _fd_grad(f, x, eps):
    g = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp[i] += eps
        xm[i] -= eps
        g[i] = (f(xp) - f(xm)) / (2 * eps)
    return g


@pytest.mark.parametrize("kind,n", [(0, 6), (1, 9), (2, 12), (3, 12), (4, 12)])
def test_fd_distance_derivatives(orc, kind, n):
    rng = np.random.default_rng(kind)
    for _ in range(5):
        x = rng.standard_normal(n)
        f = lambda y: orc.d2(kind, y)
        g, h = orc.d2_grad_hess(kind, x)
        gfd = _fd_grad(f, x, 1e-6)
        assert np.linalg.norm(g - gfd) <= 1e-6 * max(1.0, np.linalg.norm(gfd))
        hfd = np.stack([_fd_grad(lambda y: orc.d2_grad_hess(kind, y)[0][i], x, 1e-6) for i in range(n)])
        assert np.linalg.norm(h - hfd) <= 1e-5 * max(1.0, np.linalg.norm(hfd))
        assert np.allclose(h, h.T, atol=1e-12 * np.abs(h).max())


def test_fd_mollifier_reference_vertex_set(orc):
    # the vertex set and eps_x of derivTest_e (EDGE_EDGE_MOLLIFIER.h:526-580)
    x = np.array([0.0, 0.0, 0.0, 1.0, 0.1, 0.0, 0.0, 1.1, -0.1, 0.0, 0.1, -1.1])
    eps_x = 10.0
    e, g, H = orc.mollifier(x, eps_x)
    c = orc.d2(4, x)
    assert c < eps_x
    assert abs(e - (2 - c / eps_x) * c / eps_x) < 1e-15
    gfd = _fd_grad(lambda y: orc.mollifier(y, eps_x)[0], x, 1e-6)
    assert np.linalg.norm(g - gfd) <= 1e-7 * np.linalg.norm(gfd)
    hfd = np.stack([_fd_grad(lambda y: orc.mollifier(y, eps_x)[1][i], x, 1e-6) for i in range(12)])
    assert np.linalg.norm(H - hfd) <= 1e-6 * np.linalg.norm(hfd)
    # above threshold the mollifier is 1 with zero derivatives
    e1, g1, H1 = orc.mollifier(x, 1e-3)
    assert e1 == 1.0 and not g1.any() and not H1.any()


def _seg_closest_d2(p, a, b):
    ab = b - a
    t = np.clip(np.dot(p - a, ab) / np.dot(ab, ab), 0, 1)
    return np.sum((p - (a + t * ab)) ** 2)


def test_pt_type_distance_is_true_minimum(orc):
    rng = np.random.default_rng(3)
    for _ in range(400):
        x = rng.standard_normal(12)
        p, t0, t1, t2 = x.reshape(4, 3)
        dmin = orc.d2(5, x)
        # brute force: sample the triangle densely and the edges exactly
        cands = [_seg_closest_d2(p, t0, t1), _seg_closest_d2(p, t1, t2), _seg_closest_d2(p, t2, t0)]
        n = np.cross(t1 - t0, t2 - t0)
        A = np.stack([t1 - t0, t2 - t0], 1)
        uv = np.linalg.lstsq(A, p - t0, rcond=None)[0]
        if uv[0] >= 0 and uv[1] >= 0 and uv.sum() <= 1:
            cands.append(np.dot(p - t0, n) ** 2 / np.dot(n, n))
        assert abs(dmin - min(cands)) <= 1e-9 * max(1.0, min(cands))


def test_ee_type_distance_is_true_minimum(orc):
    rng = np.random.default_rng(4)
    for _ in range(400):
        x = rng.standard_normal(12)
        a0, a1, b0, b1 = x.reshape(4, 3)
        d = orc.d2(6, x)
        # dist^2 from a point of segment a to segment b is convex in the parameter:
        # ternary search gives the exact segment-segment minimum
        f = lambda s: _seg_closest_d2(a0 + s * (a1 - a0), b0, b1)
        lo, hi = 0.0, 1.0
        for _ in range(200):
            m1, m2 = lo + (hi - lo) / 3, hi - (hi - lo) / 3
            if f(m1) < f(m2):
                hi = m2
            else:
                lo = m1
        best = f(0.5 * (lo + hi))
        assert abs(d - best) <= 1e-9 * max(1.0, best)


def test_make_pd_matches_eigen_clamp(orc):
    rng = np.random.default_rng(5)
    for n in (3, 6, 9, 12):
        for _ in range(10):
            A = rng.standard_normal((n, n))
            A = A + A.T
            P = orc.make_pd(A)
            w, V = np.linalg.eigh(A)
            ref = (V * np.maximum(w, 0)) @ V.T
            assert np.abs(P - ref).max() <= 1e-10 * np.abs(A).max()
            B = A @ A.T  # PSD input: unchanged
            assert np.abs(orc.make_pd(B) - B).max() <= 1e-10 * np.abs(B).max()


def _traj_min_d2(kind, verts, disp, t_end, samples=2000):
    f = {0: 0, 1: 7, 2: 5, 3: 6}[kind]
    return min(ORC_D2(f, (verts + t * disp).ravel()) for t in np.linspace(0, t_end, samples))


def test_accd_is_conservative(orc):
    """A hit's time keeps the pair apart; a miss means no contact up to toc_in."""
    global ORC_D2
    ORC_D2 = orc.d2
    import workloads
    w = workloads.contact_pairs(400, seed=11, sep_range=(1e-3, 1e-2))
    th = 2e-4
    toc, hit, iters, ov = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], eta=0.1, thickness=th, toc_in=1.0)
    assert ov == 0
    assert hit.sum() > 0 and (hit == 0).sum() > 0
    nv = {0: 2, 1: 3, 2: 4, 3: 4}
    for i in range(0, 400, 7):
        k = int(w["type"][i])
        ids = w["idx"][i, :nv[k]]
        V, D = w["x"][ids], w["dx"][ids]
        t_end = toc[i] if hit[i] else 1.0
        assert 0 < toc[i] <= 1.0
        assert _traj_min_d2(k, V, D, t_end, 300) > th * th


def test_rod_elements_match_reference_golden(orc):
    """Rod stretching and bending derivatives (ROD_STRETCHING.h, ROD_BENDING.h) of
    the oracle's dual-number restatement against the reference's generated
    g_MS/H_MS and g_RB/H_RB on the golden inputs (unprojected Hessians)."""
    G = np.load(GOLD)
    for x, kl, g, H in zip(G["x_MS"], G["kl_MS"], G["g_MS"], G["H_MS"]):
        _, go, Ho = orc.rod_spring(x, kl[1], kl[0], project=False)
        assert np.allclose(go, g, rtol=1e-11, atol=1e-11 * np.abs(g).max())
        assert np.allclose(Ho, H, rtol=1e-10, atol=1e-10 * np.abs(H).max())
    for x, g, H in zip(G["x_RB"], G["g_RB"], G["H_RB"]):
        _, go, Ho = orc.rod_bending(x, 1.0, 1.0, project=False)
        assert np.allclose(go, g, rtol=1e-10, atol=1e-10 * np.abs(g).max())
        assert np.allclose(Ho, H, rtol=1e-9, atol=1e-9 * np.abs(H).max())

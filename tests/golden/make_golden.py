"""Generates tests/golden/reference_derivs.npz from the reference's own code.

The reference's symbolic-toolbox derivative routines (g_PT/H_PT, g_EE/H_EE,
g_PE3D/H_PE3D, g_EECN2/H_EECN2, the rod's g_MS/H_MS and g_RB/H_RB), its contact
barrier functions, its strain-limiting barrier (INEXT.h) and its friction
mollifier (FRICTION_UTILS.h), its edge-edge mollifier scalars and its
dihedral-angle derivatives are compiled from the
Codim-IPC sources by ``oracle/build.py:build_ref`` into
``oracle/_ref/libcipc_ref.so``; this script evaluates them on seeded inputs and
stores inputs and outputs, so that the oracle and the CUDA kernels can be
checked against the reference on machines without its sources.

Inputs: 48 random vertex sets per kind (standard normal coordinates) plus the
fixed vertex set of the reference's derivTest_EECross / derivTest_e
(EDGE_EDGE_MOLLIFIER.h:384-438), barrier arguments spanning 1e-12..1, and
strain-limit triples (s, limit, threshold) on both sides of 1, squared slips
on both sides of the friction mollifier's switch, 48 random hinge stencils,
32 edge pairs inside the mollifier's range and elastic-IPC barrier arguments.
Run:  python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as ob  # noqa: E402


def main():
    path = ob.build_ref()
    if path is None:
        raise SystemExit("reference sources not available")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    for n in ("ref_g_PT", "ref_H_PT", "ref_g_EE", "ref_H_EE", "ref_g_PE3D", "ref_H_PE3D", "ref_g_EECN2",
              "ref_H_EECN2"):
        getattr(L, n).argtypes = [P, P]
    L.ref_barrier.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, P]
    rng = np.random.default_rng(20210801)
    fixed = np.array([0.0, 0.0, 0.0, 1.0, 0.1, 0.0, 0.0, 1.1, -0.1, 0.0, 0.1, -1.1])
    out = {}
    for kind, n in (("PT", 12), ("EE", 12), ("PE3D", 9), ("EECN2", 12)):
        X = np.vstack([fixed[None, :], rng.standard_normal((48, 12))])
        G = np.zeros((X.shape[0], n))
        H = np.zeros((X.shape[0], n, n))
        for i, x in enumerate(X):
            xx = np.ascontiguousarray(x)
            g = np.zeros(12)
            h = np.zeros(144)
            getattr(L, "ref_g_" + kind)(xx.ctypes.data, g.ctypes.data)
            getattr(L, "ref_H_" + kind)(xx.ctypes.data, h.ctypes.data)
            G[i] = g[:n]
            H[i] = h[:n * n].reshape(n, n)
        out["x_" + kind] = X[:, :n].copy()
        out["g_" + kind] = G
        out["H_" + kind] = H
    args = []
    for d in 10.0 ** rng.uniform(-12, 0, 64):
        dhat = d * rng.uniform(1.01, 100.0)
        kappa = 10.0 ** rng.uniform(-2, 11)
        o = np.zeros(3)
        L.ref_barrier(d, dhat, kappa, o.ctypes.data)
        args.append([d, dhat, kappa, o[0], o[1], o[2]])
    out["barrier"] = np.array(args)
    # discrete rod stretching (g_MS/H_MS with E_young = k, rest length l) and
    # bending (g_RB/H_RB of |kb|^2)
    for n in ("ref_g_MS", "ref_H_MS"):
        getattr(L, n).argtypes = [ctypes.c_double, ctypes.c_double, P, P]
    for n in ("ref_g_RB", "ref_H_RB"):
        getattr(L, n).argtypes = [P, P]
    XS = rng.standard_normal((32, 6))
    KL = np.column_stack([10.0 ** rng.uniform(-1, 7, 32), rng.uniform(0.2, 2.0, 32)])
    GS = np.zeros((32, 6))
    HS = np.zeros((32, 6, 6))
    for i in range(32):
        xx = np.ascontiguousarray(XS[i])
        g = np.zeros(6)
        h = np.zeros(36)
        L.ref_g_MS(KL[i, 0], KL[i, 1], xx.ctypes.data, g.ctypes.data)
        L.ref_H_MS(KL[i, 0], KL[i, 1], xx.ctypes.data, h.ctypes.data)
        GS[i], HS[i] = g, h.reshape(6, 6)
    out.update(x_MS=XS, kl_MS=KL, g_MS=GS, H_MS=HS)
    XB = rng.standard_normal((32, 9))
    GB = np.zeros((32, 9))
    HB = np.zeros((32, 9, 9))
    for i in range(32):
        xx = np.ascontiguousarray(XB[i])
        g = np.zeros(9)
        h = np.zeros(81)
        L.ref_g_RB(xx.ctypes.data, g.ctypes.data)
        L.ref_H_RB(xx.ctypes.data, h.ctypes.data)
        GB[i], HB[i] = g, h.reshape(9, 9)
    out.update(x_RB=XB, g_RB=GB, H_RB=HB)
    # strain-limiting barrier of one singular value (INEXT.h f/g/h_sl_u for the
    # upper limit, f/g/h_sl_l for the lower), from its own seeded stream so the
    # arrays above are unchanged
    L.ref_sl.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, P]
    rs = np.random.default_rng(20240601)
    rows = []
    for _ in range(48):
        slim = 1.0 + 10.0 ** rs.uniform(-3, -0.5)
        shat = 1.0 + (slim - 1.0) * rs.uniform(0.0, 0.9)
        sv = shat + (slim - shat) * rs.uniform(0.02, 0.98)
        o = np.zeros(6)
        L.ref_sl(sv, slim, shat, o.ctypes.data)
        rows.append([0, sv, slim, shat, o[0], o[1], o[2]])
    for _ in range(48):
        slim = 1.0 - 10.0 ** rs.uniform(-3, -0.5)
        shat = 1.0 - (1.0 - slim) * rs.uniform(0.0, 0.9)
        sv = shat - (shat - slim) * rs.uniform(0.02, 0.98)
        o = np.zeros(6)
        L.ref_sl(sv, slim, shat, o.ctypes.data)
        rows.append([1, sv, slim, shat, o[3], o[4], o[5]])
    out["strain_barrier"] = np.array(rows)
    # friction mollifier (FRICTION_UTILS.h f0_SF, f1_SF_Div_RelDXNorm, f2_SF_Term)
    # on both sides of the C1 switch |u| = epsv h
    L.ref_friction.argtypes = [ctypes.c_double, ctypes.c_double, P]
    rf = np.random.default_rng(20240602)
    rows = []
    for _ in range(64):
        eh = 10.0 ** rf.uniform(-8, -2)
        x2 = (eh * 10.0 ** rf.uniform(-3, 1)) ** 2
        o = np.zeros(3)
        L.ref_friction(x2, eh, o.ctypes.data)
        rows.append([x2, eh, o[0], o[1], o[2]])
    out["friction"] = np.array(rows)
    # dihedral-angle gradient and Hessian (DIHEDRAL_ANGLE.h g_DA / H_DA, generated
    # for the unsigned acos angle) on random hinge stencils (x0, x1, x2, x3)
    L.ref_g_DA.argtypes = [P, P]
    L.ref_H_DA.argtypes = [P, P]
    rd = np.random.default_rng(20240603)
    XD = rd.standard_normal((48, 12))
    GD = np.zeros((48, 12))
    HD = np.zeros((48, 12, 12))
    for i in range(48):
        xx = np.ascontiguousarray(XD[i])
        g = np.zeros(12)
        h = np.zeros(144)
        L.ref_g_DA(xx.ctypes.data, g.ctypes.data)
        L.ref_H_DA(xx.ctypes.data, h.ctypes.data)
        GD[i], HD[i] = g, h.reshape(12, 12)
    out.update(x_DA=XD, g_DA=GD, H_DA=HD)
    # the edge-edge mollifier e(c) = EEM(c, eps_x) of c = |ea x eb|^2 with its
    # chain-rule gradient and Hessian (g_EEM / H_EEM with g_EECN2 / H_EECN2)
    L.ref_eem.argtypes = [ctypes.c_double, ctypes.c_double, P]
    rm = np.random.default_rng(20240604)
    XM = rm.standard_normal((32, 12))
    EPS = np.zeros(32)
    EM = np.zeros(32)
    GM = np.zeros((32, 12))
    HM = np.zeros((32, 12, 12))
    for i in range(32):
        xx = np.ascontiguousarray(XM[i])
        c = float(np.sum(np.cross(xx[3:6] - xx[0:3], xx[9:12] - xx[6:9]) ** 2))
        EPS[i] = c * rm.uniform(1.05, 20.0)
        o = np.zeros(3)
        L.ref_eem(c, EPS[i], o.ctypes.data)
        g = np.zeros(12)
        h = np.zeros(144)
        L.ref_g_EECN2(xx.ctypes.data, g.ctypes.data)
        L.ref_H_EECN2(xx.ctypes.data, h.ctypes.data)
        EM[i] = o[0]
        GM[i] = o[1] * g
        HM[i] = o[1] * h.reshape(12, 12) + o[2] * np.outer(g, g)
    out.update(x_EEM=XM, eps_EEM=EPS, e_EEM=EM, g_EEM=GM, H_EEM=HM)
    # the elastic-IPC branch of the barrier (Barrier<true> and its derivatives)
    L.ref_barrier_elastic.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, P]
    rb = np.random.default_rng(20240605)
    rows = []
    for d in 10.0 ** rb.uniform(-12, 0, 48):
        dhat = d * rb.uniform(1.01, 100.0)
        kappa = 10.0 ** rb.uniform(-2, 11)
        o = np.zeros(3)
        L.ref_barrier_elastic(d, dhat, kappa, o.ctypes.data)
        rows.append([d, dhat, kappa, o[0], o[1], o[2]])
    out["barrier_elastic"] = np.array(rows)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_derivs.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
